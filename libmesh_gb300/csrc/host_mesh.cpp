// Host mirror of libMesh's structured mesh generation.
//
// Produces the node coordinates, connectivity (libMesh local node order) and
// side boundary ids that a libMesh ReplicatedMesh holds after
//   MeshTools::Generation::build_cube           src/mesh/mesh_generation.C:317-1937
//   MeshTools::Modification::all_tri (HEX8)     src/mesh/mesh_modification.C:449-1180
//   MeshBase::all_second_order (TET4 -> TET10)  src/mesh/unstructured_mesh.C:60-640
// each followed by prepare_for_use(), whose ReplicatedMesh::renumber_nodes_and_elements
// (src/mesh/replicated_mesh.C:700-860) renumbers nodes in first-touch order
// over the elements.  Mesh generation is the input side of the assembly path:
// the assembly kernels never call it.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <new>

#include "lmg_internal.h"

namespace lmg {

// ------------------------------------------------------------ topology tables
// Side-to-node maps follow libMesh's ordering (src/geom/cell_hex8.C:42,
// cell_hex27.C side_nodes_map, cell_tet4.C side_nodes_map, cell_tet10.C side_nodes_map).
static const int HEX8_SIDES[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5},
                                     {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};
static const int HEX27_SIDES[6][9] = {{0, 3, 2, 1, 11, 10, 9, 8, 20},
                                      {0, 1, 5, 4, 8, 13, 16, 12, 21},
                                      {1, 2, 6, 5, 9, 14, 17, 13, 22},
                                      {2, 3, 7, 6, 10, 15, 18, 14, 23},
                                      {3, 0, 4, 7, 11, 12, 19, 15, 24},
                                      {4, 5, 6, 7, 16, 17, 18, 19, 25}};
static const int TET4_SIDES[4][3] = {{0, 2, 1}, {0, 1, 3}, {1, 2, 3}, {2, 0, 3}};
static const int TET10_SIDES[4][6] = {
    {0, 2, 1, 6, 5, 4}, {0, 1, 3, 4, 8, 7}, {1, 2, 3, 5, 9, 8}, {2, 0, 3, 6, 7, 9}};
// TET14 sides (cell_tet14.C side_nodes_map): the TET10 side and its face node.
static const int TET14_SIDES[4][7] = {
    {0, 2, 1, 6, 5, 4, 10}, {0, 1, 3, 4, 8, 7, 11}, {1, 2, 3, 5, 9, 8, 12}, {2, 0, 3, 6, 7, 9, 13}};
// PRISM6 sides (cell_prism6.C side_nodes_map): two triangles, three quads.
static const int PRISM6_SIDES[5][4] = {{0, 2, 1, -1}, {0, 1, 4, 3}, {1, 2, 5, 4}, {2, 0, 3, 5}, {3, 4, 5, -1}};
// PRISM18 / PRISM21 sides (cell_prism18.C, cell_prism21.C side_nodes_map): the
// triangles with their mid-edge nodes (and face node 18 / 19 on PRISM21), the
// quadrilaterals with mid-edge nodes and face node.
static const int PRISM21_SIDES[5][9] = {{0, 2, 1, 8, 7, 6, 18, -1, -1},
                                        {0, 1, 4, 3, 6, 10, 12, 9, 15},
                                        {1, 2, 5, 4, 7, 11, 13, 10, 16},
                                        {2, 0, 3, 5, 8, 9, 14, 11, 17},
                                        {3, 4, 5, 12, 13, 14, 19, -1, -1}};
// Vertices adjacent to TET10 mid-edge nodes 4..9 (cell_tet10.C _second_order_adjacent_vertices).
static const int TET10_EDGE_VERTS[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};

int nodes_per_elem(int t) {
  switch (t) {
    case LMG_TET4: return 4;
    case LMG_TET10: return 10;
    case LMG_TET14: return 14;
    case LMG_HEX8: return 8;
    case LMG_HEX27: return 27;
    case LMG_PRISM6: return 6;
    case LMG_PRISM18: return 18;
    case LMG_PRISM21: return 21;
    default: return 0;
  }
}
int sides_per_elem(int t) {
  switch (t) {
    case LMG_TET4: case LMG_TET10: case LMG_TET14: return 4;
    case LMG_HEX8: case LMG_HEX27: return 6;
    case LMG_PRISM6: case LMG_PRISM18: case LMG_PRISM21: return 5;
    default: return 0;
  }
}
int vertices_per_elem(int t) {
  switch (t) {
    case LMG_TET4: case LMG_TET10: case LMG_TET14: return 4;
    case LMG_HEX8: case LMG_HEX27: return 8;
    case LMG_PRISM6: case LMG_PRISM18: case LMG_PRISM21: return 6;
    default: return 0;
  }
}
int side_nodes(int t, int s, int *out) {
  switch (t) {
    case LMG_HEX8: for (int i = 0; i < 4; ++i) out[i] = HEX8_SIDES[s][i]; return 4;
    case LMG_HEX27: for (int i = 0; i < 9; ++i) out[i] = HEX27_SIDES[s][i]; return 9;
    case LMG_TET4: for (int i = 0; i < 3; ++i) out[i] = TET4_SIDES[s][i]; return 3;
    case LMG_TET10: for (int i = 0; i < 6; ++i) out[i] = TET10_SIDES[s][i]; return 6;
    case LMG_TET14: for (int i = 0; i < 7; ++i) out[i] = TET14_SIDES[s][i]; return 7;
    case LMG_PRISM6: {
      const int k = (s == 0 || s == 4) ? 3 : 4;
      for (int i = 0; i < k; ++i) out[i] = PRISM6_SIDES[s][i];
      return k;
    }
    case LMG_PRISM18:
    case LMG_PRISM21: {
      const int k = (s == 0 || s == 4) ? (t == LMG_PRISM21 ? 7 : 6) : 9;
      for (int i = 0; i < k; ++i) out[i] = PRISM21_SIDES[s][i];
      return k;
    }
    default: return 0;
  }
}

// ------------------------------------------------------------ build_cube
// Grid node index of build_cube's idx() (mesh_generation.C:118-157): a linear
// grid for HEX8, the doubled grid for HEX27.
static inline int64_t grid_idx(int64_t gx, int64_t gy, int64_t i, int64_t j, int64_t k) {
  return i + gx * (j + k * gy);
}

// PRISM6 build_cube (mesh_generation.C:1501-1545): the HEX8 node grid, two
// prisms per grid cell split along the (i+1, j) - (i, j+1) diagonal, in
// k, j, i cell order; side ids on the triangles (0 bottom, 5 top) and on the
// quads that lie on the cube faces.
static std::string build_cube_prism6(HostMesh &m, int nx, int ny, int nz) {
  const int64_t gx = (int64_t)nx + 1, gy = (int64_t)ny + 1, gz = (int64_t)nz + 1;
  m.elem_type = LMG_PRISM6;
  m.npe = 6;
  m.nsides = 5;
  m.xyz.resize((size_t)(gx * gy * gz) * 3);
  for (int64_t k = 0; k < gz; ++k)
    for (int64_t j = 0; j < gy; ++j)
      for (int64_t i = 0; i < gx; ++i) {
        const int64_t id = grid_idx(gx, gy, i, j, k);
        m.xyz[3 * id + 0] = (double)i / (double)nx * (1.0 - 0.0) + 0.0;
        m.xyz[3 * id + 1] = (double)j / (double)ny * (1.0 - 0.0) + 0.0;
        m.xyz[3 * id + 2] = (double)k / (double)nz * (1.0 - 0.0) + 0.0;
      }
  const int64_t E = 2 * (int64_t)nx * ny * nz;
  m.conn.resize((size_t)(E * 6));
  m.side_bid.assign((size_t)(E * 5), (int8_t)-1);
  int64_t e = 0;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        int32_t *c = &m.conn[(size_t)(e * 6)];
        int8_t *sb = &m.side_bid[(size_t)(e * 5)];
        c[0] = (int32_t)grid_idx(gx, gy, i, j, k);
        c[1] = (int32_t)grid_idx(gx, gy, i + 1, j, k);
        c[2] = (int32_t)grid_idx(gx, gy, i, j + 1, k);
        c[3] = (int32_t)grid_idx(gx, gy, i, j, k + 1);
        c[4] = (int32_t)grid_idx(gx, gy, i + 1, j, k + 1);
        c[5] = (int32_t)grid_idx(gx, gy, i, j + 1, k + 1);
        if (i == 0) sb[3] = 4;
        if (j == 0) sb[1] = 1;
        if (k == 0) sb[0] = 0;
        if (k == nz - 1) sb[4] = 5;
        ++e;
        c = &m.conn[(size_t)(e * 6)];
        sb = &m.side_bid[(size_t)(e * 5)];
        c[0] = (int32_t)grid_idx(gx, gy, i + 1, j, k);
        c[1] = (int32_t)grid_idx(gx, gy, i + 1, j + 1, k);
        c[2] = (int32_t)grid_idx(gx, gy, i, j + 1, k);
        c[3] = (int32_t)grid_idx(gx, gy, i + 1, j, k + 1);
        c[4] = (int32_t)grid_idx(gx, gy, i + 1, j + 1, k + 1);
        c[5] = (int32_t)grid_idx(gx, gy, i, j + 1, k + 1);
        if (i == nx - 1) sb[1] = 2;
        if (j == ny - 1) sb[2] = 3;
        if (k == 0) sb[0] = 0;
        if (k == nz - 1) sb[4] = 5;
        ++e;
      }
  renumber_nodes_first_touch(m);
  return "";
}

// PRISM18 / PRISM21 build_cube (mesh_generation.C:1324-1377, 1634-1745): the
// doubled node grid, for PRISM21 followed by two triangle-centre nodes per grid
// cell on each of the 2 nz + 1 levels, at ((i + 1/3) / nx, (j + 1/3) / ny) and
// ((i + 2/3) / nx, (j + 2/3) / ny); two prisms per cell as for PRISM6, with
// their mid-edge nodes, quad-face nodes and (PRISM21) triangle-face and
// interior nodes taken from the grid.
static std::string build_cube_prism_hi(HostMesh &m, int nx, int ny, int nz, int type) {
  const int64_t gx = 2 * (int64_t)nx + 1, gy = 2 * (int64_t)ny + 1, gz = 2 * (int64_t)nz + 1;
  const bool p21 = type == LMG_PRISM21;
  const int npe = p21 ? 21 : 18;
  m.elem_type = type;
  m.npe = npe;
  m.nsides = 5;
  const int64_t n_grid = gx * gy * gz, n_tri = p21 ? gz * (int64_t)nx * ny * 2 : 0;
  m.xyz.resize((size_t)(n_grid + n_tri) * 3);
  for (int64_t k = 0; k < gz; ++k)
    for (int64_t j = 0; j < gy; ++j)
      for (int64_t i = 0; i < gx; ++i) {
        const int64_t id = grid_idx(gx, gy, i, j, k);
        m.xyz[3 * id + 0] = (double)i / (double)(2 * nx) * (1.0 - 0.0) + 0.0;
        m.xyz[3 * id + 1] = (double)j / (double)(2 * ny) * (1.0 - 0.0) + 0.0;
        m.xyz[3 * id + 2] = (double)k / (double)(2 * nz) * (1.0 - 0.0) + 0.0;
      }
  if (p21) {
    const double kmax = (double)(2 * nz);
    int64_t id = n_grid;
    for (int64_t k = 0; k < gz; ++k)
      for (int64_t j = 0; j < ny; ++j)
        for (int64_t i = 0; i < nx; ++i)
          for (int t = 1; t <= 2; ++t, ++id) {
            const double third = (double)t / 3.0;
            m.xyz[3 * id + 0] = ((double)i + third) / (double)nx * (1.0 - 0.0) + 0.0;
            m.xyz[3 * id + 1] = ((double)j + third) / (double)ny * (1.0 - 0.0) + 0.0;
            m.xyz[3 * id + 2] = (double)k / kmax * (1.0 - 0.0) + 0.0;
          }
  }
  const int64_t E = 2 * (int64_t)nx * ny * nz;
  m.conn.resize((size_t)(E * npe));
  m.side_bid.assign((size_t)(E * 5), (int8_t)-1);
  // grid offsets (i, j, k) of nodes 0..17 of the first and second prism of a cell
  static const int A[18][3] = {{0, 0, 0}, {2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {2, 0, 2}, {0, 2, 2},
                               {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 1}, {0, 2, 1},
                               {1, 0, 2}, {1, 1, 2}, {0, 1, 2}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
  static const int B[18][3] = {{2, 0, 0}, {2, 2, 0}, {0, 2, 0}, {2, 0, 2}, {2, 2, 2}, {0, 2, 2},
                               {2, 1, 0}, {1, 2, 0}, {1, 1, 0}, {2, 0, 1}, {2, 2, 1}, {0, 2, 1},
                               {2, 1, 2}, {1, 2, 2}, {1, 1, 2}, {2, 1, 1}, {1, 2, 1}, {1, 1, 1}};
  int64_t e = 0;
  for (int k = 0; k < 2 * nz; k += 2)
    for (int j = 0; j < 2 * ny; j += 2)
      for (int i = 0; i < 2 * nx; i += 2)
        for (int second = 0; second < 2; ++second, ++e) {
          const int (*off)[3] = second ? B : A;
          int32_t *c = &m.conn[(size_t)(e * npe)];
          for (int a = 0; a < 18; ++a) c[a] = (int32_t)grid_idx(gx, gy, i + off[a][0], j + off[a][1], k + off[a][2]);
          if (p21) {  // triangle-face nodes 18 (bottom), 19 (top) and interior node 20
            const int64_t cell = (int64_t)(j / 2) * nx + i / 2;
            c[18] = (int32_t)(n_grid + ((int64_t)k * nx * ny + cell) * 2 + second);
            c[19] = (int32_t)(n_grid + ((int64_t)(k + 2) * nx * ny + cell) * 2 + second);
            c[20] = (int32_t)(n_grid + ((int64_t)(k + 1) * nx * ny + cell) * 2 + second);
          }
          int8_t *sb = &m.side_bid[(size_t)(e * 5)];
          if (!second) {
            if (i == 0) sb[3] = 4;
            if (j == 0) sb[1] = 1;
          } else {
            if (i == 2 * (nx - 1)) sb[1] = 2;
            if (j == 2 * (ny - 1)) sb[2] = 3;
          }
          if (k == 0) sb[0] = 0;
          if (k == 2 * (nz - 1)) sb[4] = 5;
        }
  renumber_nodes_first_touch(m);
  return "";
}

std::string build_cube_hex(HostMesh &m, int nx, int ny, int nz, int type) {
  if (nx <= 0 || ny <= 0 || nz <= 0) return "build_cube: nx, ny, nz must be positive";
  if (type != LMG_HEX8 && type != LMG_HEX27 && type != LMG_PRISM6 && type != LMG_PRISM18 && type != LMG_PRISM21)
    return "build_cube: type must be HEX8, HEX27, PRISM6, PRISM18 or PRISM21";
  if (type == LMG_PRISM6) return build_cube_prism6(m, nx, ny, nz);
  if (type == LMG_PRISM18 || type == LMG_PRISM21) return build_cube_prism_hi(m, nx, ny, nz, type);
  const int f = (type == LMG_HEX8) ? 1 : 2;  // grid refinement factor
  const int64_t gx = (int64_t)f * nx + 1, gy = (int64_t)f * ny + 1, gz = (int64_t)f * nz + 1;
  m.elem_type = type;
  m.npe = nodes_per_elem(type);
  m.nsides = 6;
  m.xyz.resize((size_t)(gx * gy * gz) * 3);
  // Nodes in k, j, i loop order; coordinate = (i / (f*nx)) * (xmax - xmin) + xmin
  // with the unit cube, i.e. exactly i / (f*nx) (mesh_generation.C:1281-1377, 1776-1786).
  for (int64_t k = 0; k < gz; ++k)
    for (int64_t j = 0; j < gy; ++j)
      for (int64_t i = 0; i < gx; ++i) {
        const int64_t id = grid_idx(gx, gy, i, j, k);
        double x = (double)i / (double)(f * nx);
        double y = (double)j / (double)(f * ny);
        double z = (double)k / (double)(f * nz);
        m.xyz[3 * id + 0] = x * (1.0 - 0.0) + 0.0;
        m.xyz[3 * id + 1] = y * (1.0 - 0.0) + 0.0;
        m.xyz[3 * id + 2] = z * (1.0 - 0.0) + 0.0;
      }
  const int64_t E = (int64_t)nx * ny * nz;
  m.conn.resize((size_t)(E * m.npe));
  m.side_bid.assign((size_t)(E * 6), (int8_t)-1);
  int64_t e = 0;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i, ++e) {
        int32_t *c = &m.conn[(size_t)(e * m.npe)];
        if (type == LMG_HEX8) {
          // mesh_generation.C:1398-1430
          c[0] = (int32_t)grid_idx(gx, gy, i, j, k);
          c[1] = (int32_t)grid_idx(gx, gy, i + 1, j, k);
          c[2] = (int32_t)grid_idx(gx, gy, i + 1, j + 1, k);
          c[3] = (int32_t)grid_idx(gx, gy, i, j + 1, k);
          c[4] = (int32_t)grid_idx(gx, gy, i, j, k + 1);
          c[5] = (int32_t)grid_idx(gx, gy, i + 1, j, k + 1);
          c[6] = (int32_t)grid_idx(gx, gy, i + 1, j + 1, k + 1);
          c[7] = (int32_t)grid_idx(gx, gy, i, j + 1, k + 1);
        } else {
          // HEX27 on the doubled grid, mesh_generation.C:1569-1604
          const int I = 2 * i, J = 2 * j, K = 2 * k;
          static const int off[27][3] = {
              {0, 0, 0}, {2, 0, 0}, {2, 2, 0}, {0, 2, 0}, {0, 0, 2}, {2, 0, 2}, {2, 2, 2},
              {0, 2, 2}, {1, 0, 0}, {2, 1, 0}, {1, 2, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 1},
              {2, 2, 1}, {0, 2, 1}, {1, 0, 2}, {2, 1, 2}, {1, 2, 2}, {0, 1, 2}, {1, 1, 0},
              {1, 0, 1}, {2, 1, 1}, {1, 2, 1}, {0, 1, 1}, {1, 1, 2}, {1, 1, 1}};
          for (int a = 0; a < 27; ++a)
            c[a] = (int32_t)grid_idx(gx, gy, I + off[a][0], J + off[a][1], K + off[a][2]);
        }
        int8_t *sb = &m.side_bid[(size_t)(e * 6)];
        if (k == 0) sb[0] = 0;
        if (k == nz - 1) sb[5] = 5;
        if (j == 0) sb[1] = 1;
        if (j == ny - 1) sb[3] = 3;
        if (i == 0) sb[4] = 4;
        if (i == nx - 1) sb[2] = 2;
      }
  renumber_nodes_first_touch(m);
  return "";
}

// ReplicatedMesh::renumber_nodes_and_elements (replicated_mesh.C:700-860):
// nodes receive ids in order of first appearance over elements (in element id
// order, local node order); untouched nodes keep their relative order after.
void renumber_nodes_first_touch(HostMesh &m) {
  const int64_t N = m.n_nodes();
  std::vector<int32_t> newid((size_t)N, -1);
  int32_t next = 0;
  for (size_t p = 0; p < m.conn.size(); ++p) {
    int32_t &slot = newid[(size_t)m.conn[p]];
    if (slot < 0) slot = next++;
  }
  for (int64_t n = 0; n < N; ++n)
    if (newid[(size_t)n] < 0) newid[(size_t)n] = next++;
  std::vector<double> xyz((size_t)N * 3);
  for (int64_t n = 0; n < N; ++n)
    for (int d = 0; d < 3; ++d) xyz[(size_t)(3 * newid[(size_t)n] + d)] = m.xyz[(size_t)(3 * n + d)];
  m.xyz.swap(xyz);
  for (auto &c : m.conn) c = newid[(size_t)c];
}

// Interior vertices of a unit-cube grid move by U[-amp*h, amp*h] per
// coordinate, in node id order, three draws per interior node.
void jitter_interior(HostMesh &m, double amp, int nx, int ny, int nz, uint64_t seed) {
  if (amp == 0.0) return;
  SplitMix64 rng(seed);
  const double h[3] = {1.0 / nx, 1.0 / ny, 1.0 / nz};
  const int64_t N = m.n_nodes();
  for (int64_t n = 0; n < N; ++n) {
    double *p = &m.xyz[(size_t)(3 * n)];
    bool interior = true;
    for (int d = 0; d < 3; ++d)
      if (p[d] == 0.0 || p[d] == 1.0) interior = false;
    if (!interior) continue;
    for (int d = 0; d < 3; ++d) p[d] += (2.0 * rng.u01() - 1.0) * amp * h[d];
  }
}

}  // namespace lmg
