// Reference-element tables for the element kernels: QGauss points and weights,
// LAGRANGE shape values and reference gradients at those points, and the
// reference tensors used by the affine fast path.  Built once per
// (element type, FE order, quadrature order) on the host and uploaded.
//
// Rules follow libMesh's QGauss (src/quadrature/quadrature_gauss_1D.C:30-80,
// src/quadrature/quadrature_gauss_3D.C:30-226, src/quadrature/quadrature.C:283-305):
// an order-p rule integrates degree-p polynomials exactly, hexes use the
// tensor product with the first coordinate fastest, tets use the published
// Zienkiewicz-Taylor (orders 1-3) and Keast (order 4, 11 points, one negative
// weight) rules.  The 1D Gauss-Legendre nodes are computed here by Newton
// iteration on P_n in long double.
#include <cmath>

#include "lmg_internal.h"

namespace lmg {

namespace {

void gauss_legendre(int np, std::vector<double> &x, std::vector<double> &w) {
  x.assign(np, 0.0);
  w.assign(np, 0.0);
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int i = 0; i < np; ++i) {
    // i-th node from the left: cos(pi (np - i - 0.25) / (np + 0.5)) start.
    long double z = cosl(pi * (np - i - 0.25L) / (np + 0.5L));
    long double dp = 0;
    for (int it = 0; it < 100; ++it) {
      long double p0 = 1, p1 = z;
      for (int k = 2; k <= np; ++k) {
        long double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      if (np == 1) { p1 = z; p0 = 1; }
      dp = np * (z * p1 - p0) / (z * z - 1);
      long double dz = p1 / dp;
      z -= dz;
      if (fabsl(dz) < 1e-30L) break;
    }
    long double p0 = 1, p1 = z;
    for (int k = 2; k <= np; ++k) {
      long double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    dp = (np == 1) ? 1.0L : np * (z * p1 - p0) / (z * z - 1);
    x[i] = (double)z;
    w[i] = (double)(2.0L / ((1 - z * z) * dp * dp));
  }
  // 3-5 points: the 32-digit values libMesh tabulates (quadrature_gauss_1D.C:30-120),
  // so that difference quotients taken at these points match bit for bit.
  if (np == 3) {
    x[0] = -7.7459666924148337703585307995648e-01;
    w[0] = 5.0 / 9;
    w[1] = 8.0 / 9;
  } else if (np == 4) {
    x[0] = -8.6113631159405257522394648889281e-01;
    x[1] = -3.3998104358485626480266575910324e-01;
    w[0] = 3.4785484513745385737306394922200e-01;
    w[1] = 6.5214515486254614262693605077800e-01;
  } else if (np == 5) {
    x[0] = -9.0617984593866399279762687829939e-01;
    x[1] = -5.3846931010568309103631442070021e-01;
    w[0] = 2.3692688505618908751426404071992e-01;
    w[1] = 4.7862867049936646804129151483564e-01;
    w[2] = 5.6888888888888888888888888888889e-01;
  }
  if (np % 2 == 1) x[np / 2] = 0.0;  // the middle node is exactly zero
  for (int i = 0; i < np / 2; ++i) {  // exact symmetry, as libMesh stores it
    x[np - 1 - i] = -x[i];
    w[np - 1 - i] = w[i];
  }
}

void tet_rule(int order, std::vector<double> &p, std::vector<double> &w) {
  p.clear();
  w.clear();
  auto add = [&](double a, double b, double c, double wt) {
    p.push_back(a); p.push_back(b); p.push_back(c); w.push_back(wt);
  };
  if (order <= 1) {
    add(0.25, 0.25, 0.25, 1.0 / 6.0);
  } else if (order == 2) {
    const double b = 0.25 * (1.0 - std::sqrt(5.0) / 5.0), a = 1.0 - 3.0 * b;
    add(a, b, b, 1.0 / 24); add(b, a, b, 1.0 / 24); add(b, b, a, 1.0 / 24); add(b, b, b, 1.0 / 24);
  } else if (order == 3) {
    add(0.25, 0.25, 0.25, -2.0 / 15.0);
    add(0.5, 1.0 / 6, 1.0 / 6, 0.075); add(1.0 / 6, 0.5, 1.0 / 6, 0.075);
    add(1.0 / 6, 1.0 / 6, 0.5, 0.075); add(1.0 / 6, 1.0 / 6, 1.0 / 6, 0.075);
  } else if (order == 5) {
    // Walkington's 14-point degree-5 rule (quadrature_gauss_3D.C:231-287): two
    // 4-orbits (a, a, a), (a, b, a), (b, a, a), (a, a, b) with b = 1 - 3a, and
    // a 6-orbit with b = (1 - 2a) / 2, in the reference's point order.
    const double a[3] = {0.31088591926330060980, 0.092735250310891226402, 0.045503704125649649492};
    const double wt[3] = {0.018781320953002641800, 0.012248840519393658257, 0.0070910034628469110730};
    for (int i = 0; i < 2; ++i) {
      const double b = 1. - 3. * a[i];
      add(a[i], a[i], a[i], wt[i]); add(a[i], b, a[i], wt[i]); add(b, a[i], a[i], wt[i]); add(a[i], a[i], b, wt[i]);
    }
    const double b = 0.5 * (1. - 2. * a[2]), c = a[2], w6 = wt[2];
    add(b, b, c, w6); add(b, c, c, w6); add(c, c, b, w6); add(c, b, c, w6); add(b, c, b, w6); add(c, b, b, w6);
  } else if (order == 6) {
    // Keast's 24-point degree-6 rule (quadrature_gauss_3D.C:401-420 through
    // keast_rule, quadrature_gauss.C:43-180): three 4-orbits (a, b, b),
    // (b, a, b), (b, b, a), (b, b, b) and one 12-orbit, with the reference's
    // 18-digit values.
    const double r[3][3] = {{0.356191386222544953e+00, 0.214602871259151684e+00, 0.00665379170969464506e+00},
                            {0.877978124396165982e+00, 0.0406739585346113397e+00, 0.00167953517588677620e+00},
                            {0.0329863295731730594e+00, 0.322337890142275646e+00, 0.00922619692394239843e+00}};
    for (int i = 0; i < 3; ++i) {
      const double a = r[i][0], b = r[i][1], wt = r[i][2];
      add(a, b, b, wt); add(b, a, b, wt); add(b, b, a, wt); add(b, b, b, wt);
    }
    const double a = 0.0636610018750175299e+00, b = 0.269672331458315867e+00, c = 0.603005664791649076e+00,
                 wt = 0.00803571428571428248e+00;
    add(a, a, b, wt); add(a, a, c, wt); add(b, a, a, wt); add(c, a, a, wt); add(a, b, a, wt); add(a, c, a, wt);
    add(a, b, c, wt); add(a, c, b, wt); add(b, a, c, wt); add(b, c, a, wt); add(c, a, b, wt); add(c, b, a, wt);
  } else if (order == 4) {
    // Keast (1986) degree-4 rule: centroid, a 4-orbit and a 6-orbit, with the
    // 18-digit values libMesh tabulates (quadrature_gauss_3D.C:198-226), so
    // that difference quotients of shapes at these points agree bit for bit.
    add(0.25, 0.25, 0.25, -0.131555555555555556e-01);
    const double a4 = 0.785714285714285714e+00, b4 = 0.714285714285714285e-01, w4 = 0.762222222222222222e-02;
    add(a4, b4, b4, w4); add(b4, a4, b4, w4); add(b4, b4, a4, w4); add(b4, b4, b4, w4);
    const double a6 = 0.399403576166799219e+00, b6 = 0.100596423833200785e+00, w6 = 0.248888888888888889e-01;
    add(a6, a6, b6, w6); add(a6, b6, b6, w6); add(b6, b6, a6, w6);
    add(b6, a6, b6, w6); add(b6, a6, a6, w6); add(a6, b6, a6, w6);
  }
}

// Triangle QGauss rules on the reference triangle (0,0), (1,0), (0,1), as
// libMesh tabulates them (src/quadrature/quadrature_gauss_2D.C:73-260): the
// centroid (FIRST), the three interior points (SECOND), the 4-point conical
// product rule (THIRD), the published Dunavant rule of degree 4 (6 points) and
// the degree-5 rule (7 points), expanded from their orbits in the same point
// order.  The
// literal values are kept so that a point's difference quotients agree bit for
// bit with the reference's.
void tri_rule(int order, std::vector<double> &p, std::vector<double> &w) {
  p.clear();
  w.clear();
  auto add = [&](double a, double b, double wt) { p.push_back(a); p.push_back(b); w.push_back(wt); };
  // Dunavant orbit expansion: a 1-orbit at the centroid, a 3-orbit (a, a, 1-2a)
  // in the order (a, a), (a, 1-2a), (1-2a, a).
  auto orbit = [&](double a, double wt) {
    add(a, a, wt);
    add(a, 1.0 - 2.0 * a, wt);
    add(1.0 - 2.0 * a, a, wt);
  };
  if (order <= 1) {
    add(1.0 / 3, 1.0 / 3, 0.5);
  } else if (order == 2) {
    add(2.0 / 3, 1.0 / 6, 1.0 / 6); add(1.0 / 6, 2.0 / 3, 1.0 / 6); add(1.0 / 6, 1.0 / 6, 1.0 / 6);
  } else if (order == 3) {
    add(1.5505102572168219018027159252941e-01, 1.7855872826361642311703513337422e-01, 1.5902069087198858469718450103758e-01);
    add(6.4494897427831780981972840747059e-01, 7.5031110222608118177475598324603e-02, 9.0979309128011415302815498962418e-02);
    add(1.5505102572168219018027159252941e-01, 6.6639024601470138670269327409637e-01, 1.5902069087198858469718450103758e-01);
    add(6.4494897427831780981972840747059e-01, 2.8001991549907407200279599420481e-01, 9.0979309128011415302815498962418e-02);
  } else if (order == 4) {
    orbit(4.4594849091596488631832925388305e-01, 1.1169079483900573284750350421656e-01);
    orbit(9.1576213509770743459571463402202e-02, 5.4975871827660933819163162450105e-02);
  } else {  // degree 5 (Walkington): centroid and two 3-orbits given in closed form
    add(1.0 / 3, 1.0 / 3, 9.0 / 80);
    orbit(2.0 / 7 + std::sqrt(15.0) / 21, 31.0 / 480 + std::sqrt(15.0) / 2400);
    orbit(2.0 / 7 - std::sqrt(15.0) / 21, 31.0 / 480 - std::sqrt(15.0) / 2400);
  }
}

// Hex node -> 1D index tables (the node numbering of libMesh's HEX8 / HEX27).
const int HEX8_I[3][8] = {{0, 1, 1, 0, 0, 1, 1, 0}, {0, 0, 1, 1, 0, 0, 1, 1}, {0, 0, 0, 0, 1, 1, 1, 1}};
const int HEX27_I[3][27] = {
    {0, 1, 1, 0, 0, 1, 1, 0, 2, 1, 2, 0, 0, 1, 1, 0, 2, 1, 2, 0, 2, 2, 1, 2, 0, 2, 2},
    {0, 0, 1, 1, 0, 0, 1, 1, 0, 2, 1, 2, 0, 0, 1, 1, 0, 2, 1, 2, 2, 0, 2, 1, 2, 2, 2},
    {0, 0, 0, 0, 1, 1, 1, 1, 0, 0, 0, 0, 2, 2, 2, 2, 1, 1, 1, 1, 0, 2, 2, 2, 2, 1, 2}};

void l1d(int order, int i, double x, double &v, double &d) {
  if (order == 1) {
    v = (i == 0) ? 0.5 * (1.0 - x) : 0.5 * (1.0 + x);
    d = (i == 0) ? -0.5 : 0.5;
  } else {
    if (i == 0) { v = 0.5 * x * (x - 1.0); d = x - 0.5; }
    else if (i == 1) { v = 0.5 * x * (x + 1.0); d = x + 0.5; }
    else { v = 1.0 - x * x; d = -2.0 * x; }
  }
}

// Values and reference gradients of the n LAGRANGE shapes at point p.
int lagrange_shapes(int type, int order, const double *p, double *v, double *g) {
  if (type == LMG_HEX8 || type == LMG_HEX27) {
    const int n = (order == 1) ? 8 : 27;
    if (order == 2 && type != LMG_HEX27) return 0;
    for (int a = 0; a < n; ++a) {
      double s[3], ds[3];
      for (int m = 0; m < 3; ++m) {
        const int idx = (order == 1) ? HEX8_I[m][a] : HEX27_I[m][a];
        l1d(order, idx, p[m], s[m], ds[m]);
      }
      v[a] = s[0] * s[1] * s[2];
      g[3 * a + 0] = ds[0] * s[1] * s[2];
      g[3 * a + 1] = s[0] * ds[1] * s[2];
      g[3 * a + 2] = s[0] * s[1] * ds[2];
    }
    return n;
  }
  if (type == LMG_PRISM6) {
    // fe_lagrange_shape_3D.C PRISM6: TRI3 shape (1 - xi - eta, xi, eta) times
    // the 1-D linear shape in zeta; nodes 0-2 at zeta = -1, 3-5 at zeta = +1.
    if (order != 1) return 0;
    const double t[3] = {1. - p[0] - p[1], p[0], p[1]};
    const double dt[3][2] = {{-1., -1.}, {1., 0.}, {0., 1.}};
    for (int a = 0; a < 6; ++a) {
      const int i1 = a % 3, i0 = a / 3;
      const double l = i0 == 0 ? .5 * (1. - p[2]) : .5 * (1. + p[2]), dl = i0 == 0 ? -.5 : .5;
      v[a] = t[i1] * l;
      g[3 * a + 0] = dt[i1][0] * l;
      g[3 * a + 1] = dt[i1][1] * l;
      g[3 * a + 2] = t[i1] * dl;
    }
    return 6;
  }
  if (type == LMG_TET4 || type == LMG_TET10 || type == LMG_TET14) {
    const double z[4] = {1.0 - p[0] - p[1] - p[2], p[0], p[1], p[2]};
    const double dz[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    if (order == 1) {
      for (int a = 0; a < 4; ++a) {
        v[a] = z[a];
        for (int m = 0; m < 3; ++m) g[3 * a + m] = dz[a][m];
      }
      return 4;
    }
    if (type == LMG_TET14) {
      // TET14 (fe_lagrange_shape_3D.C:1402-1460, derivatives :2931-3260):
      // quadratic functions corrected by the face bubbles z_a z_b z_c.
      const double b[4] = {z[0] * z[1] * z[2], z[0] * z[1] * z[3], z[1] * z[2] * z[3], z[0] * z[2] * z[3]};
      // d bubble / d xi_j for bubbles 012, 013, 123, 023
      const double db[3][4] = {{(z[0] - z[1]) * z[2], (z[0] - z[1]) * z[3], z[2] * z[3], -z[2] * z[3]},
                               {(z[0] - z[2]) * z[1], -z[1] * z[3], z[1] * z[3], (z[0] - z[2]) * z[3]},
                               {-z[1] * z[2], (z[0] - z[3]) * z[1], z[1] * z[2], (z[0] - z[3]) * z[2]}};
      static const int VB[4][3] = {{0, 1, 3}, {0, 1, 2}, {0, 3, 2}, {1, 3, 2}};  // bubbles at each vertex
      static const int EN[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
      static const int EB[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 3}, {1, 2}, {3, 2}};  // bubbles at each edge
      static const int FB[4] = {0, 1, 2, 3};
      for (int a = 0; a < 4; ++a) {
        v[a] = z[a] * (2. * z[a] - 1.) + 3. * (b[VB[a][0]] + b[VB[a][1]] + b[VB[a][2]]);
        for (int m = 0; m < 3; ++m)
          g[3 * a + m] = (4. * z[a] - 1.) * dz[a][m] + 3. * (db[m][VB[a][0]] + db[m][VB[a][1]] + db[m][VB[a][2]]);
      }
      for (int k = 0; k < 6; ++k) {
        const int i = EN[k][0], j = EN[k][1];
        // node 6 is written 4 z2 z0 in the reference
        v[4 + k] = (k == 2 ? 4. * z[2] * z[0] : 4. * z[i] * z[j]) - 12. * (b[EB[k][0]] + b[EB[k][1]]);
        for (int m = 0; m < 3; ++m)
          g[3 * (4 + k) + m] = 4. * (z[i] * dz[j][m] + dz[i][m] * z[j]) - 12. * (db[m][EB[k][0]] + db[m][EB[k][1]]);
      }
      for (int f = 0; f < 4; ++f) {
        v[10 + f] = 27. * b[FB[f]];
        for (int m = 0; m < 3; ++m) g[3 * (10 + f) + m] = 27. * db[m][FB[f]];
      }
      return 14;
    }
    if (type != LMG_TET10) return 0;
    static const int EV[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
    for (int a = 0; a < 4; ++a) {
      v[a] = z[a] * (2.0 * z[a] - 1.0);
      for (int m = 0; m < 3; ++m) g[3 * a + m] = (4.0 * z[a] - 1.0) * dz[a][m];
    }
    for (int k = 0; k < 6; ++k) {
      const int i = EV[k][0], j = EV[k][1];
      v[4 + k] = 4.0 * z[i] * z[j];
      for (int m = 0; m < 3; ++m) g[3 * (4 + k) + m] = 4.0 * (z[i] * dz[j][m] + dz[i][m] * z[j]);
    }
    return 10;
  }
  return 0;
}

// fe_hierarchic_1D_shape (src/fe/fe_hierarchic_shape_1D.C:430-498): linear
// end functions, then (xi^i - 1)/i! (even i) and (xi^i - xi)/i! (odd i).
double hier1d(int i, double xi) {
  switch (i) {
    case 0: return .5 * (1. - xi);
    case 1: return .5 * (1. + xi);
    case 2: return (xi * xi - 1.) / 2.;
    default: return (xi * xi * xi - xi) / 6.;
  }
}

// HIERARCHIC hex shapes for p <= 2 (fe_hierarchic_shape_3D.C:2249-2290 with
// cube_indices, :166-760): the tensor index of dof i is the HEX27 node index
// table (vertices, one edge dof per edge, one dof per face, one interior dof).
// The bases are even in every coordinate, so the reflections of cube_indices
// leave them unchanged, but its face swaps move coordinates between the
// product's factors: at SECOND order the shapes follow the element's
// orientation pattern (hex27_p2_shape, given its vertices X8).  Value = (s0 s1) s2;
// derivative = (shape(p + eps e_j) - shape(p - eps e_j)) / 2. / eps with
// eps = 1e-6 (fe_fdm_deriv, src/fe/fe.C:794-811, 929-944).
//
// Tets (TET4 FIRST, TET10 SECOND): barycentric vertex functions and, per edge
// (v0, v1) of the TET4 edge list, c^2 * hier1d(2, (z1 - z0) / c) with
// c = z0 + z1 ((z1 - z0)^2 / 2 where c is exactly 0); std::pow as the
// reference evaluates it, so the difference quotients match bit for bit.
double hier_tet(int a, const double *x) {
  const double zeta[4] = {1 - x[0] - x[1] - x[2], x[0], x[1], x[2]};
  if (a < 4) return zeta[a];
  static const int EN[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
  const unsigned k = 2;
  const double c = zeta[EN[a - 4][0]] + zeta[EN[a - 4][1]], num = zeta[EN[a - 4][1]] - zeta[EN[a - 4][0]];
  if (c == 0.) return std::pow(num, k) / 2u;
  const double flip = 1;
  return flip * std::pow(c, k) * hier1d(2, num / c);
}

//
// PRISM6 FIRST (prism_indices vertices): TRI vertex function times the 1-D
// end function, the same products as LAGRANGE; derivatives by the same
// difference quotient.
double hier_prism6(int a, const double *x) {
  const double t[3] = {1. - x[0] - x[1], x[0], x[1]};
  const int i01 = a % 3, i2 = a / 3;
  return t[i01] * (i2 == 0 ? .5 * (1. - x[2]) : .5 * (1. + x[2]));
}

int hierarchic_shapes(int type, int order, const double *p, double *v, double *g, const double *X8) {
  const bool tet = (type == LMG_TET4 && order == 1) || (type == LMG_TET10 && order == 2);
  const bool tet3 = false;  // cubic tets depend on the element: hier_tet3_shapes
  const bool prism = type == LMG_PRISM6 && order == 1;
  if (!((type == LMG_HEX8 && order == 1) || (type == LMG_HEX27 && order == 2) || tet || prism) || tet3) return 0;
  const int n = prism ? 6 : tet ? (order == 1 ? 4 : 10) : (order == 1) ? 8 : 27;
  auto shape = [&](int a, const double *x) {
    if (prism) return hier_prism6(a, x);
    if (tet) return hier_tet(a, x);
    if (order == 2 && X8) return hex27_p2_shape(reinterpret_cast<const double(*)[3]>(X8), a, x);
    const int i0 = (order == 1) ? HEX8_I[0][a] : HEX27_I[0][a], i1 = (order == 1) ? HEX8_I[1][a] : HEX27_I[1][a],
              i2 = (order == 1) ? HEX8_I[2][a] : HEX27_I[2][a];
    return hier1d(i0, x[0]) * hier1d(i1, x[1]) * hier1d(i2, x[2]);
  };
  const double eps = 1.e-6;
  for (int a = 0; a < n; ++a) {
    v[a] = shape(a, p);
    for (int j = 0; j < 3; ++j) {
      double pp[3] = {p[0], p[1], p[2]}, pm[3] = {p[0], p[1], p[2]};
      pp[j] += eps;
      pm[j] -= eps;
      g[3 * a + j] = (shape(a, pp) - shape(a, pm)) / 2. / eps;
    }
  }
  return n;
}

}  // namespace

// Cubic HIERARCHIC tets (FEType{THIRD, HIERARCHIC} on TET14,
// fe_hierarchic_shape_3D.C:2361-2440): vertices; per edge e the bases of
// order 2 and 3, c^order * hier1d(order, (z1 - z0) / c) with c = z0 + z1
// ((z1 - z0)^order / order! where c is exactly 0), the order-3 one negated
// when positive_edge_orientation(e) holds (elem.C:3634-3640: the edge's first
// vertex is lexicographically greater); per face f the bubble
// ((1 * z_a) * z_b) * z_c over the face's vertices as orient_triangle sorts
// them (fe_hierarchic_shape_3D.C:2193-2243).
TetOrient tet_orient(const double *X) {
  auto greater = [&](int a, int b) {  // TypeVector::operator> (type_vector.C:95-105)
    for (int d = 0; d < 3; ++d) {
      if (X[3 * a + d] > X[3 * b + d]) return true;
      if (X[3 * a + d] < X[3 * b + d]) return false;
    }
    return false;
  };
  static const int EN[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
  static const int SV[4][3] = {{0, 2, 1}, {0, 1, 3}, {1, 2, 3}, {2, 0, 3}};  // Tet4 side vertices
  TetOrient o;
  o.flip = 0;
  for (int e = 0; e < 6; ++e)
    if (greater(EN[e][0], EN[e][1])) o.flip |= (uint8_t)(1u << e);
  for (int f = 0; f < 4; ++f) {
    int v[3] = {SV[f][0], SV[f][1], SV[f][2]};
    bool lastcheck = true;
    if (greater(v[0], v[1])) { std::swap(v[0], v[1]); lastcheck = true; }
    if (greater(v[1], v[2])) std::swap(v[1], v[2]);
    if (lastcheck && greater(v[0], v[1])) std::swap(v[0], v[1]);
    for (int k = 0; k < 3; ++k) o.fv[f][k] = (uint8_t)v[k];
  }
  return o;
}

static double hier_tet3(const TetOrient &o, int a, const double *x) {
  const double zeta[4] = {1 - x[0] - x[1] - x[2], x[0], x[1], x[2]};
  if (a < 4) return zeta[a];
  static const int EN[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
  if (a < 16) {
    const int edge = (a - 4) / 2;
    const unsigned basisorder = (unsigned)(a - 2 - 2 * edge);
    double flip = 1;
    if (basisorder % 2 && ((o.flip >> edge) & 1u)) flip = -1;
    const double c = zeta[EN[edge][0]] + zeta[EN[edge][1]], num = zeta[EN[edge][1]] - zeta[EN[edge][0]];
    if (c == 0.) {
      unsigned fact = 1;
      for (unsigned n = 2; n <= basisorder; ++n) fact *= n;
      return std::pow(num, basisorder) / fact;
    }
    return flip * std::pow(c, basisorder) * hier1d((int)basisorder, num / c);
  }
  const int f = a - 16;
  double r = 1;
  r *= zeta[o.fv[f][0]];
  r *= zeta[o.fv[f][1]];
  r *= zeta[o.fv[f][2]];
  return r;
}

int hier_tet3_shapes(const TetOrient &o, const double *p, double *v, double *g) {
  const double eps = 1.e-6;
  for (int a = 0; a < 20; ++a) {
    v[a] = hier_tet3(o, a, p);
    for (int j = 0; j < 3; ++j) {
      double pp[3] = {p[0], p[1], p[2]}, pm[3] = {p[0], p[1], p[2]};
      pp[j] += eps;
      pm[j] -= eps;
      g[3 * a + j] = (hier_tet3(o, a, pp) - hier_tet3(o, a, pm)) / 2. / eps;
    }
  }
  return 20;
}

std::string build_fe_tables(FETables &t, int type, int fe_order, int q_order, int family, const double *X8) {
  t = FETables();
  t.elem_type = type;
  t.fe_order = fe_order;
  t.q_order = q_order;
  t.family = family;
  if (fe_order < 1 || fe_order > 2) return "fe_order must be FIRST or SECOND";
  if (family != 0 && family != 1) return "unknown FE family";
  if (family == 1 && !((type == LMG_HEX8 && fe_order == 1) || (type == LMG_HEX27 && fe_order == 2) ||
                       (type == LMG_TET4 && fe_order == 1) || (type == LMG_TET10 && fe_order == 2) ||
                       (type == LMG_PRISM6 && fe_order == 1)))
    return "HIERARCHIC is built for FIRST on HEX8 / TET4 / PRISM6 and SECOND on HEX27 / TET10";
  auto fe_shapes = [&](const double *p, double *v, double *g) {
    return family == 1 ? hierarchic_shapes(type, fe_order, p, v, g, X8) : lagrange_shapes(type, fe_order, p, v, g);
  };
  const bool hex = (type == LMG_HEX8 || type == LMG_HEX27);
  const bool tet = (type == LMG_TET4 || type == LMG_TET10 || type == LMG_TET14);
  const bool prism = type == LMG_PRISM6;
  if (!hex && !tet && !prism) return "unsupported element type";
  const int geo_order = (type == LMG_HEX27 || type == LMG_TET10) ? 2 : type == LMG_TET14 ? 3 : 1;
  if (hex) {
    std::vector<double> x, w;
    gauss_legendre(q_order / 2 + 1, x, w);
    const int np = (int)x.size();
    for (int k = 0; k < np; ++k)
      for (int j = 0; j < np; ++j)
        for (int i = 0; i < np; ++i) {
          t.qp.push_back(x[i]); t.qp.push_back(x[j]); t.qp.push_back(x[k]);
          t.qw.push_back(w[i] * w[j] * w[k]);
        }
  } else if (prism) {
    // tensor_product_prism (quadrature.C:310-331): triangle point fastest,
    // then the 1-D Gauss point in zeta.
    if (q_order > 5) return "prism quadrature above FIFTH is not built";
    std::vector<double> x, w, tp, tw;
    gauss_legendre(q_order / 2 + 1, x, w);
    tri_rule(q_order, tp, tw);
    for (size_t j = 0; j < x.size(); ++j)
      for (size_t i = 0; i < tw.size(); ++i) {
        t.qp.push_back(tp[2 * i]); t.qp.push_back(tp[2 * i + 1]); t.qp.push_back(x[j]);
        t.qw.push_back(tw[i] * w[j]);
      }
  } else {
    if (q_order > 6) return "tet quadrature above SIXTH is not built";
    tet_rule(q_order, t.qp, t.qw);
  }
  t.q = (int)t.qw.size();
  double v[27], g[81];
  t.n = fe_shapes(&t.qp[0], v, g);
  t.n_geo = lagrange_shapes(type, geo_order, &t.qp[0], v, g);
  if (!t.n || !t.n_geo) return "unsupported element type / order";
  t.phi.resize((size_t)t.q * t.n);
  t.dphi.resize((size_t)t.q * t.n * 3);
  t.gphi.resize((size_t)t.q * t.n_geo);
  t.gdphi.resize((size_t)t.q * t.n_geo * 3);
  for (int q = 0; q < t.q; ++q) {
    fe_shapes(&t.qp[3 * q], v, g);
    for (int a = 0; a < t.n; ++a) {
      t.phi[(size_t)q * t.n + a] = v[a];
      for (int m = 0; m < 3; ++m) t.dphi[((size_t)q * t.n + a) * 3 + m] = g[3 * a + m];
    }
    lagrange_shapes(type, geo_order, &t.qp[3 * q], v, g);
    for (int a = 0; a < t.n_geo; ++a) {
      t.gphi[(size_t)q * t.n_geo + a] = v[a];
      for (int m = 0; m < 3; ++m) t.gdphi[((size_t)q * t.n_geo + a) * 3 + m] = g[3 * a + m];
    }
  }
  const int n = t.n;
  t.S.assign((size_t)9 * n * n, 0.0);
  t.M.assign((size_t)n * n, 0.0);
  for (int q = 0; q < t.q; ++q)
    for (int a = 0; a < n; ++a)
      for (int b = 0; b < n; ++b) {
        t.M[(size_t)a * n + b] += t.qw[q] * t.phi[(size_t)q * n + a] * t.phi[(size_t)q * n + b];
        for (int m = 0; m < 3; ++m)
          for (int mm = 0; mm < 3; ++mm)
            t.S[(((size_t)(m * 3 + mm) * n) + a) * n + b] +=
                t.qw[q] * t.dphi[((size_t)q * n + a) * 3 + m] * t.dphi[((size_t)q * n + b) * 3 + mm];
      }
  return "";
}

namespace {
// libMesh relative_fuzzy_equals on 3-vectors (include/utils/fuzzy_equals.h:78-84):
// l1(a - b) <= tol * (l1(a) + l1(b)), with affine_tol = TOLERANCE^2 = 1e-12.
bool rfe_tol(const double *a, const double *b, double tol) {
  double d = 0, na = 0, nb = 0;
  for (int i = 0; i < 3; ++i) {
    d += std::fabs(a[i] - b[i]);
    na += std::fabs(a[i]);
    nb += std::fabs(b[i]);
  }
  return d <= tol * (na + nb);
}
bool rfe(const double *a, const double *b) {
  const double tol = 1e-6 * 1e-6;
  double d = 0, na = 0, nb = 0;
  for (int i = 0; i < 3; ++i) {
    d += std::fabs(a[i] - b[i]);
    na += std::fabs(a[i]);
    nb += std::fabs(b[i]);
  }
  return d <= tol * (na + nb);
}
void sub(const double *P, int i, int j, double *o) {
  for (int d = 0; d < 3; ++d) o[d] = P[3 * i + d] - P[3 * j + d];
}
}  // namespace

bool elem_has_affine_map(int type, const double *P) {
  double v[3], w[3];
  switch (type) {
    case LMG_PRISM6: {  // cell_prism6.C:199-207: the three z edges are parallel translates
      sub(P, 3, 0, v);
      sub(P, 4, 1, w); if (!rfe(v, w)) return false;
      sub(P, 5, 2, w); return rfe(v, w);
    }
    case LMG_PRISM18:    // cell_prism18.C:122-150
    case LMG_PRISM21: {  // cell_prism21.C:139-180: straight edges, then centred triangle-face nodes
      sub(P, 3, 0, v);
      sub(P, 4, 1, w); if (!rfe(v, w)) return false;
      sub(P, 5, 2, w); if (!rfe(v, w)) return false;
      for (int d = 0; d < 3; ++d) v[d] /= 2;
      static const int Z[6][2] = {{9, 0}, {10, 1}, {11, 2}, {15, 6}, {16, 7}, {17, 8}};
      for (auto &z : Z) {
        sub(P, z[0], z[1], w);
        if (!rfe(v, w)) return false;
      }
      static const int T[3][4] = {{1, 0, 6, 0}, {2, 0, 8, 0}, {2, 1, 7, 1}};  // v = (b - a) / 2 against m - a, m' - a'
      for (auto &t : T) {
        sub(P, t[0], t[1], v);
        for (int d = 0; d < 3; ++d) v[d] /= 2;
        sub(P, t[2], t[3], w); if (!rfe(v, w)) return false;
        sub(P, t[2] + 6, t[3] + 3, w); if (!rfe(v, w)) return false;
      }
      if (type == LMG_PRISM18) return true;
      static const int F[3][4] = {{2, 1, 0, 18}, {5, 4, 3, 19}, {11, 10, 9, 20}};  // c + b - 2 a against 3 (m - a)
      for (auto &f : F) {
        for (int d = 0; d < 3; ++d) {
          v[d] = P[3 * f[0] + d] + P[3 * f[1] + d] - 2 * P[3 * f[2] + d];
          w[d] = (P[3 * f[3] + d] - P[3 * f[2] + d]) * 3;
        }
        if (!rfe_tol(v, w, 1e-6)) return false;
      }
      return true;
    }
    case LMG_TET4:
      return true;
    case LMG_TET10:    // cell_tet10.C:143-172
    case LMG_TET14: {  // cell_tet14.C:153-194: straight edges, then midface nodes
      static const int E[6][3] = {{1, 0, 4}, {2, 1, 5}, {2, 0, 6}, {3, 0, 7}, {3, 1, 8}, {3, 2, 9}};
      for (int k = 0; k < 6; ++k) {
        sub(P, E[k][0], E[k][1], v);
        sub(P, E[k][2], E[k][1], w);
        for (int d = 0; d < 3; ++d) w[d] *= 2;
        if (!rfe(v, w)) return false;
      }
      if (type == LMG_TET10) return true;
      // (v_b0 + v_c0) against 3 (p_face - p_0), with v_ij = p_i - p_j
      static const int F[4][5] = {{2, 0, 1, 0, 10}, {3, 0, 1, 0, 11}, {3, 1, 2, 1, 12}, {3, 0, 2, 0, 13}};
      double a[3], b[3];
      for (int f = 0; f < 4; ++f) {
        sub(P, F[f][0], F[f][1], a);
        sub(P, F[f][2], F[f][3], b);
        const int base = f == 2 ? 1 : 0;
        for (int d = 0; d < 3; ++d) v[d] = a[d] + b[d];
        sub(P, F[f][4], base, w);
        for (int d = 0; d < 3; ++d) w[d] *= 3;
        if (!rfe(v, w)) return false;
      }
      return true;
    }
    case LMG_HEX8: {  // cell_hex8.C:121-135
      sub(P, 1, 0, v);
      sub(P, 2, 3, w); if (!rfe(v, w)) return false;
      sub(P, 5, 4, w); if (!rfe(v, w)) return false;
      sub(P, 6, 7, w); if (!rfe(v, w)) return false;
      sub(P, 4, 0, v);
      sub(P, 7, 3, w); return rfe(v, w);
    }
    case LMG_HEX27: {  // cell_hex27.C:125-170
      sub(P, 1, 0, v);
      sub(P, 2, 3, w); if (!rfe(v, w)) return false;
      sub(P, 5, 4, w); if (!rfe(v, w)) return false;
      sub(P, 6, 7, w); if (!rfe(v, w)) return false;
      for (int d = 0; d < 3; ++d) v[d] /= 2;
      static const int X[9][2] = {{8, 0}, {10, 3}, {16, 4}, {18, 7}, {20, 11},
                                  {21, 12}, {23, 15}, {25, 19}, {26, 24}};
      for (auto &p : X) { sub(P, p[0], p[1], w); if (!rfe(v, w)) return false; }
      sub(P, 4, 0, v);
      sub(P, 7, 3, w); if (!rfe(v, w)) return false;
      for (int d = 0; d < 3; ++d) v[d] /= 2;
      static const int Z[6][2] = {{12, 0}, {13, 1}, {14, 2}, {15, 3}, {22, 9}, {24, 11}};
      for (auto &p : Z) { sub(P, p[0], p[1], w); if (!rfe(v, w)) return false; }
      sub(P, 3, 0, v);
      for (int d = 0; d < 3; ++d) v[d] /= 2;
      static const int Y[4][2] = {{11, 0}, {9, 1}, {17, 5}, {19, 4}};
      for (auto &p : Y) { sub(P, p[0], p[1], w); if (!rfe(v, w)) return false; }
      return true;
    }
    default:
      return false;
  }
}

}  // namespace lmg
