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
// Refinement tree of a structured hex cube (host_amr.cpp).  Every element
// ever created keeps its id (children are appended, as MeshRefinement::add_elem
// does); node and element corners live on an integer lattice whose level-0
// element edge is AMR_S0, so coincident nodes are found exactly.
constexpr int64_t AMR_S0 = 1024;
constexpr int AMR_MAX_LEVEL = 8;
struct AmrTree {
  bool on = false;
  int nx = 0, ny = 0, nz = 0;
  std::vector<int32_t> conn;          // [n_all][npe], current node ids
  std::vector<int32_t> parent;        // -1 on level 0
  std::vector<int32_t> first_child;   // -1 while active
  std::vector<int8_t> level;
  std::vector<int64_t> origin;        // [n_all][3] lattice position of vertex 0
  std::vector<int8_t> side_bid;       // [n_all][6]
  std::vector<int64_t> node_lat;      // [n_nodes][3]
  std::vector<int32_t> active;        // active element ids, id order
  int64_t n_all() const { return (int64_t)parent.size(); }
};

struct HostMesh {
  int elem_type = 0;
  int npe = 0;           // nodes per element
  int nsides = 0;        // sides per element
  std::vector<double> xyz;      // [n_nodes][3]
  std::vector<int32_t> conn;    // [n_elem][npe]
  std::vector<int8_t> side_bid; // [n_elem][nsides], -1 = interior
  int cube[3] = {0, 0, 0};      // build_cube grid of an unjittered hex cube (else 0)
  AmrTree amr;                  // refinement tree once lmg_mesh_refine ran
  int64_t n_nodes() const { return (int64_t)xyz.size() / 3; }
  int64_t n_elem() const { return npe ? (int64_t)conn.size() / npe : 0; }
};

// Builders (host_mesh.cpp).  Each returns an error string, empty on success.
std::string build_cube_hex(HostMesh &m, int nx, int ny, int nz, int type);
void renumber_nodes_first_touch(HostMesh &m);
void jitter_interior(HostMesh &m, double amp, int nx, int ny, int nz, uint64_t seed);
std::string all_tri_hex8(HostMesh &m);
std::string all_second_order_tet4(HostMesh &m);

// AMR (host_amr.cpp).  amr_refine runs `cycles` rounds of: flag
// floor(fraction * n_active) random active elements, enforce the level-one
// rule across faces, refine; HostMesh::conn / side_bid then hold the active
// elements in id order.
std::string amr_refine(HostMesh &m, int cycles, double fraction, uint64_t seed);
// Constraint rows of the dofs of hanging nodes (lagrange_compute_constraints)
// for LAGRANGE variables on the active mesh, then empty rows for the dofs in
// `dirichlet` that are still free, then chain expansion (process_constraints).
// rows: dof -> (dof -> coefficient), both ascending.
struct ConstraintRows {
  std::vector<int32_t> dofs;                 // constrained dofs, ascending
  std::vector<int64_t> ptr;                  // [dofs.size() + 1]
  std::vector<int32_t> col;
  std::vector<double> val;
};
std::string amr_constraint_rows(const HostMesh &m, int n_vars, const int32_t *elem_dofs, int64_t n_dofs,
                                const uint8_t *dirichlet, ConstraintRows &out);
// The hanging-node rows formed on the device (amr_rows.cu): dof d's row has
// cnt[d] entries (-1: none) at col / val[d * width ..]; the Dirichlet rows,
// process_constraints and the output follow on the host as above.
std::string constraint_rows_from_raw(int64_t n_dofs, const int32_t *cnt, const int32_t *col, const double *val,
                                     int width, const uint8_t *dirichlet, ConstraintRows &out);
std::string amr_raw_rows_device(const HostMesh &m, int device, int n_vars, const int32_t *elem_dofs, int64_t n_dofs,
                                std::vector<int32_t> &cnt, std::vector<int32_t> &col, std::vector<double> &val);
constexpr int AMR_ROW_WIDTH = 9;  // entries of a raw hanging-node row (QUAD9 side)
// distribute_dofs on the device (dofs_device.cu): the numbering and dof_indices
// of lmg_dofmap_distribute_fe; returns an error message or "".
std::string distribute_dofs_device(int device, int64_t n_nodes, int64_t n_elem, int elem_type, const int32_t *conn,
                                   int n_vars, int fe_order, int64_t &n_dofs, int32_t *elem_dofs);

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
  int family = 0;  // 0 LAGRANGE, 1 HIERARCHIC
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
// family 1 (HIERARCHIC, hexahedra, p <= 2): products of the 1-D hierarchic
// shapes, reference derivatives by libMesh's central differences (eps = 1e-6).
// X8: for HIERARCHIC SECOND on HEX27, the vertex coordinates [8][3] of an
// element whose orientation pattern every element of the mesh shares (the
// tables then follow that pattern's evaluation order).
std::string build_fe_tables(FETables &t, int elem_type, int fe_order, int q_order, int family = 0,
                            const double *X8 = nullptr);

// Cubic HIERARCHIC hex tables (hier3_tables.cpp): each element's 64 shape
// variants and the tables over the variants that occur.
struct Hier3Tables {
  int N = 64, G = 27;            // dofs and map nodes per element
  int V = 0;                     // variants
  int q = 0;                     // quadrature points
  std::vector<uint16_t> var;     // [n_elem][64] variant of each shape
  std::vector<double> D;         // [V][V][6] affine reference tensors
  std::vector<double> M;         // [V][27]   sum_q w phi_v phi^geo_g
  std::vector<double> gd0;       // [27][3]   HEX27 map derivatives at qp 0
  // Elements grouped by their 64-variant pattern: per pattern the tensors in
  // the element's own shape order, the elements sorted by pattern, and
  // batches of at most 8 elements of one pattern.
  int P = 0;
  std::vector<double> Dp;        // [P][6][N*N]
  std::vector<double> Mp;        // [P][N][G]
  std::vector<int32_t> order;    // [n_elem] element ids sorted by pattern (stable)
  std::vector<int32_t> batch;    // [n_batch][3]: pattern, first index in order, count
};
std::string build_hier3_tables(Hier3Tables &h, int q_order, int64_t n_elem, const double *xyz, const int32_t *conn);
// HIERARCHIC SECOND on HEX27 (cube_indices at totalorder 2): the orientation
// pattern of an element from its vertex coordinates, and shape a at p as the
// reference evaluates it on such an element.
uint64_t hex27_p2_pattern(const double (*X)[3]);
double hex27_p2_shape(const double (*X)[3], int a, const double *p);

// Orientation of a TET14 for the cubic HIERARCHIC basis: bit e of flip set
// when edge e's order-3 basis is negated, fv[f] the vertices of face f as
// orient_triangle sorts them.
struct TetOrient {
  uint8_t flip = 0;
  uint8_t fv[4][3] = {};
  uint32_t key() const {
    uint32_t k = flip;
    for (int f = 0; f < 4; ++f) k = (k << 6) | (uint32_t)(fv[f][0] << 4) | (uint32_t)(fv[f][1] << 2) | fv[f][2];
    return k;
  }
};
TetOrient tet_orient(const double *X /* [4][3] vertex coordinates */);
// values [20] and reference gradients [20][3] (central differences, eps = 1e-6)
int hier_tet3_shapes(const TetOrient &o, const double *p, double *v, double *g);
std::string build_tet3_tables(Hier3Tables &h, int q_order, int64_t n_elem, const double *xyz, const int32_t *conn);
// HIERARCHIC of order 2 on PRISM18 or 3 on PRISM21 (npe = 18 / 21 nodes per
// connectivity row): the same tables over the elements' orientation records,
// with the six vertices' PRISM6 basis for the map and the load.
std::string build_prism_tables(Hier3Tables &h, int order, int q_order, int64_t n_elem, const double *xyz,
                               const int32_t *conn, int npe);

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
// Sparsity of a constrained system (DofMap::compute_sparsity with
// find_connected_dofs): every element couples the sorted union of its dofs and,
// transitively, the dofs that constrain them.  cons_ptr [n_dofs+1] / cons_col
// give each dof's constraint row (empty for free and Dirichlet dofs).
void build_constrained_graph(int64_t n_elem, int nl, const int32_t *elem_dofs, int64_t n_dofs,
                             const int64_t *cons_ptr, const int32_t *cons_col,
                             std::vector<int64_t> &row_ptr, std::vector<int32_t> &cols, int n_threads);
void build_block_graph(int64_t n_elem, int nb_per_elem, const int32_t *elem_blocks,
                       int64_t n_blocks, std::vector<int64_t> &row_ptr,
                       std::vector<int32_t> &cols, int n_threads);

}  // namespace lmg

// The opaque mesh handle of the C ABI.
struct lmg_mesh {
  lmg::HostMesh m;
  // constraint rows of the last lmg_constraint_rows call and its input checksum
  lmg::ConstraintRows rows;
  uint64_t rows_key = 0;
  bool rows_valid = false;
};
