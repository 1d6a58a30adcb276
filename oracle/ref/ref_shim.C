// Test infrastructure (oracle/_ref): the few definitions the compiled
// reference sources need from files that cannot be compiled here (libmesh.C
// and elem.C pull in the parallel library, whose submodule is absent).
// Restated from those files; every other unresolved symbol is a stub that
// aborts with its name when called (generated by oracle/ref_build.py).
#include "libmesh/elem.h"

#include <iostream>

namespace libMesh {

// libmesh.C: the library's output streams.
OStreamProxy out(std::cout);
OStreamProxy err(std::cerr);

// elem.C, Elem::positive_edge_orientation: an edge is positive when the point
// of its first node compares greater than that of its second.
bool Elem::positive_edge_orientation(const unsigned int i) const {
  return this->point(this->local_edge_node(i, 0)) > this->point(this->local_edge_node(i, 1));
}

// elem.C, Elem::positive_face_orientation: around the face's smallest vertex
// (by point comparison), the face is positive when the previous vertex
// compares less than the next one.  N, the face's vertex count, is 3 for
// triangular sides (3, 6 or 7 nodes) and 4 for quadrilateral ones.
bool Elem::positive_face_orientation(const unsigned int i) const {
  const std::vector<unsigned int> nodes = this->nodes_on_side(i);
  const unsigned int N = (nodes.size() == 3 || nodes.size() == 6 || nodes.size() == 7) ? 3 : 4;
  auto less = [&](unsigned int m, unsigned int n) { return this->point(m) < this->point(n); };
  unsigned int v = 0;
  for (unsigned int k = 1; k < N; ++k)
    if (less(nodes[k], nodes[v])) v = k;
  return less(nodes[(v + N - 1) % N], nodes[(v + 1) % N]);
}

// elem.C, Elem::set_interior_parent: the interior parent link sits after the
// element's side-neighbor links.
void Elem::set_interior_parent(Elem *p) { _elemlinks[1 + this->n_sides()] = p; }

}  // namespace libMesh
