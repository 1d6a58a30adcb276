// Internal declarations shared by the host (C++) and device (CUDA) parts of
// libmesh_gb300.  Not part of the C ABI.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/libmesh_gb300.h"

namespace lmg {

// ---------------------------------------------------------------- topology
int nodes_per_elem(int elem_type);   // 0 if unknown
int sides_per_elem(int elem_type);
int vertices_per_elem(int elem_type);
// Local node numbers on side s of elem_type (libMesh side_nodes_map order);
// returns the count written to out (out must hold 9).
int side_nodes(int elem_type, int s, int *out);

// ---------------------------------------------------------------- mesh
struct HostMesh {
  int elem_type = 0;
  int npe = 0;           // nodes per element
  int nsides = 0;        // sides per element
  std::vector<double> xyz;      // [n_nodes][3]
  std::vector<int32_t> conn;    // [n_elem][npe]
  std::vector<int8_t> side_bid; // [n_elem][nsides], -1 = interior
  int64_t n_nodes() const { return (int64_t)xyz.size() / 3; }
  int64_t n_elem() const { return npe ? (int64_t)conn.size() / npe : 0; }
};

// Builders (host_mesh.cpp).  Each returns an error string, empty on success.
std::string build_cube_hex(HostMesh &m, int nx, int ny, int nz, int type);
void renumber_nodes_first_touch(HostMesh &m);
void jitter_interior(HostMesh &m, double amp, int nx, int ny, int nz, uint64_t seed);
std::string all_tri_hex8(HostMesh &m);
std::string all_second_order_tet4(HostMesh &m);

// ---------------------------------------------------------------- rng
// splitmix64; u01 maps the top 53 bits to [0,1).
struct SplitMix64 {
  uint64_t s;
  explicit SplitMix64(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double u01() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// ---------------------------------------------------------------- FE tables
// Reference-element data for one (element type, FE order, quadrature order).
struct FETables {
  int elem_type = 0, fe_order = 0, q_order = 0;
  int n = 0;       // shape functions
  int q = 0;       // quadrature points
  int n_geo = 0;   // mapping shape functions (element default order)
  std::vector<double> qp;        // [q][3]
  std::vector<double> qw;        // [q]
  std::vector<double> phi;       // [q][n]
  std::vector<double> dphi;      // [q][n][3]  d phi / d xi_m
  std::vector<double> gphi;      // [q][n_geo]  mapping shape values
  std::vector<double> gdphi;     // [q][n_geo][3] mapping shape derivatives
  std::vector<double> S;         // [3][3][n][n]: sum_q w dphi_a/dxi_m dphi_b/dxi_n
  std::vector<double> M;         // [n][n]: sum_q w phi_a phi_b
};
std::string build_fe_tables(FETables &t, int elem_type, int fe_order, int q_order);

// libMesh Elem::has_affine_map for one element (cell_hex8.C:121, cell_hex27.C:125,
// cell_tet4 always, cell_tet10.C:143).
bool elem_has_affine_map(int elem_type, const double *pts /* [npe][3] */);

// ---------------------------------------------------------------- sparsity
// Block graph of the element-dof coupling: elements couple every block they
// touch (block = dof / bs).  row_ptr has n_blocks+1 entries, cols sorted.
// Detects node-interleaved variables (dof = bs*block + var for every element
// node) and fills elem_blocks [n_elem][nb]; bs = n_vars and nb = npe when the
// layout holds, else bs = 1 and nb = n_vars*npe (every dof is a block).
void block_structure(int64_t n_elem, int npe, int n_vars, const int32_t *elem_dofs, int &bs, int &nb,
                     std::vector<int32_t> &elem_blocks);
void build_block_graph(int64_t n_elem, int nb_per_elem, const int32_t *elem_blocks,
                       int64_t n_blocks, std::vector<int64_t> &row_ptr,
                       std::vector<int32_t> &cols, int n_threads);

}  // namespace lmg
