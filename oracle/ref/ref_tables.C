// Test infrastructure (oracle/_ref): evaluates the reference's own QGauss
// rules and LAGRANGE / HIERARCHIC shape functions.  Commands on standard
// input, results on standard output (%.17g, exact for doubles):
//   qgauss TYPE ORDER                      -> n, then n lines "x y z w"
//   lagrange TYPE ORDER N NP  p_1..p_NP    -> phi[i][q] (N*NP), dphi[c][i][q] (3*N*NP)
//   hierarchic TYPE ORDER N NN x_1..x_NN NP p_1..p_NP
//                                          -> the same for FE<3,HIERARCHIC> on an
//                                             element of TYPE with node points x
// TYPE and ORDER are libMesh's ElemType and Order values.
#include "libmesh/cell_hex27.h"
#include "libmesh/cell_hex8.h"
#include "libmesh/cell_prism18.h"
#include "libmesh/cell_prism20.h"
#include "libmesh/cell_prism21.h"
#include "libmesh/cell_prism6.h"
#include "libmesh/cell_tet10.h"
#include "libmesh/cell_tet14.h"
#include "libmesh/cell_tet4.h"
#include "libmesh/fe.h"
#include "libmesh/node.h"
#include "libmesh/quadrature_gauss.h"

#include <cstdio>
#include <iostream>
#include <memory>
#include <string>
#include <vector>

using namespace libMesh;

namespace {

std::unique_ptr<Elem> make_elem(ElemType t) {
  switch (t) {
    case HEX8: return std::make_unique<Hex8>();
    case HEX27: return std::make_unique<Hex27>();
    case TET4: return std::make_unique<Tet4>();
    case TET10: return std::make_unique<Tet10>();
    case TET14: return std::make_unique<Tet14>();
    case PRISM6: return std::make_unique<Prism6>();
    case PRISM18: return std::make_unique<Prism18>();
    case PRISM20: return std::make_unique<Prism20>();
    case PRISM21: return std::make_unique<Prism21>();
    default: return nullptr;
  }
}

std::vector<Point> read_points(int n) {
  std::vector<Point> p((size_t)n);
  for (auto &x : p) std::cin >> x(0) >> x(1) >> x(2);
  return p;
}

}  // namespace

int main() {
  std::string cmd;
  while (std::cin >> cmd) {
    int type = 0, order = 0;
    std::cin >> type >> order;
    const ElemType t = static_cast<ElemType>(type);
    const Order o = static_cast<Order>(order);
    if (cmd == "qgauss") {
      QGauss q(3, o);
      q.init(t, 0, true);
      std::printf("%u\n", q.n_points());
      for (unsigned int i = 0; i < q.n_points(); ++i)
        std::printf("%.17g %.17g %.17g %.17g\n", q.qp(i)(0), q.qp(i)(1), q.qp(i)(2), q.w(i));
    } else if (cmd == "lagrange" || cmd == "hierarchic") {
      int n = 0;
      std::cin >> n;
      std::unique_ptr<Elem> el;
      std::vector<std::unique_ptr<Node>> nodes;
      if (cmd == "hierarchic") {
        int nn = 0;
        std::cin >> nn;
        el = make_elem(t);
        if (!el || (int)el->n_nodes() != nn) {
          std::printf("error\n");
          return 1;
        }
        const std::vector<Point> X = read_points(nn);
        for (int a = 0; a < nn; ++a) {
          nodes.emplace_back(new Node(X[(size_t)a], (dof_id_type)a));
          el->set_node(a, nodes.back().get());
        }
      }
      int np = 0;
      std::cin >> np;
      const std::vector<Point> P = read_points(np);
      for (int i = 0; i < n; ++i)
        for (int q = 0; q < np; ++q)
          std::printf("%.17g\n", el ? FE<3, HIERARCHIC>::shape(el.get(), o, i, P[(size_t)q], true)
                                    : FE<3, LAGRANGE>::shape(t, o, i, P[(size_t)q]));
      for (int c = 0; c < 3; ++c)
        for (int i = 0; i < n; ++i)
          for (int q = 0; q < np; ++q)
            std::printf("%.17g\n", el ? FE<3, HIERARCHIC>::shape_deriv(el.get(), o, i, c, P[(size_t)q], true)
                                      : FE<3, LAGRANGE>::shape_deriv(t, o, i, c, P[(size_t)q]));
    } else {
      std::printf("error\n");
      return 1;
    }
    std::fflush(stdout);
  }
  return 0;
}
