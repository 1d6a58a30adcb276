// Hanging-node constraint rows on the device (lagrange_compute_constraints,
// src/fe/fe_lagrange.C:867-1063, for h-refined structured hex cubes).
//
// libMesh visits, per variable, every active element with a parent and every
// side of that child that lies on the parent's side and faces a coarser
// neighbour; each node of the child's side whose dof is not one of the parent
// side's dofs gets the row  u_node = sum_j phi_j(xi, eta) u_{parent side node j}
// (phi the parent side's LAGRANGE shapes, entries kept when
// 1e-5 < |phi| < 0.999), the first visit of a dof writing its row.  Here one
// thread takes one (variable, active element, side):
//   k_node_dofs  dof of every (node, variable) from the active elements' dof lists;
//   k_visits<false>  every candidate (dof, visit) claims its dof with atomicMin
//                on the visit's position in libMesh's loop order, so the first
//                visit wins whatever the thread schedule;
//   k_visits<true>   the winning visits write their rows (the side shapes at the
//                node's parent-side coordinates, exact lattice ratios), each
//                in ascending column order.
// The tree queries (the active element across a side) descend the refinement
// tree from the level-0 cell by lattice position, as the host's locate does.
// The arithmetic is unfused (__dmul_rn, __dadd_rn) in the host's order, so the
// rows are the host's bit for bit; the Dirichlet rows and process_constraints
// (dof_map_constraints.C:4341-4490, a sequential substitution over the few
// rows that refer to constrained dofs) follow on the host.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "lmg_internal.h"

namespace lmg {

namespace {

struct TreeArgs {
  int nx, ny, nz, npe, n_vars, ns;
  int64_t n_active, n_dofs;
  const int32_t *tconn;       // [n_all][npe] all elements' nodes
  const int32_t *parent, *first_child;
  const int8_t *level;
  const int64_t *origin;      // [n_all][3]
  const int64_t *node_lat;    // [n_nodes][3]
  const int32_t *active;      // [n_active] tree ids of the active elements
  const int32_t *node_dof;    // [n_nodes][n_vars]
  unsigned long long *claim;  // [n_dofs] first visit of each dof
  int32_t *cnt;               // [n_dofs] row length (-1: no row)
  int32_t *col;               // [n_dofs][AMR_ROW_WIDTH]
  double *val;
  int *status;
};

__constant__ int c_sides[6][9];    // side node maps of the element type (HEX8: 4, HEX27: 9)
__constant__ int c_hex8[6][4];     // HEX8 side vertices (children on a side)
__constant__ int c_vbits[8][3];    // hex vertex offsets
__constant__ int c_axis[6], c_sign[6];

__device__ int32_t d_locate(const TreeArgs &t, const int64_t p[3]) {
  const int64_t n[3] = {t.nx, t.ny, t.nz};
  int64_t c[3];
  for (int d = 0; d < 3; ++d) {
    if (p[d] <= 0 || p[d] >= n[d] * AMR_S0) return -1;
    c[d] = p[d] / AMR_S0;
  }
  int32_t e = (int32_t)(c[0] + t.nx * (c[1] + t.ny * c[2]));
  for (int depth = 0; depth < 60 && t.first_child[e] >= 0; ++depth) {
    const int64_t h = (AMR_S0 >> t.level[e]) / 2;
    int b[3];
    for (int d = 0; d < 3; ++d) b[d] = (p[d] - t.origin[3 * (int64_t)e + d]) >= h ? 1 : 0;
    int child = 0;
    for (int v = 0; v < 8; ++v)
      if (c_vbits[v][0] == b[0] && c_vbits[v][1] == b[1] && c_vbits[v][2] == b[2]) child = v;
    e = t.first_child[e] + child;
  }
  return e;
}

__device__ int32_t d_across(const TreeArgs &t, int32_t e, int s) {
  const int64_t S = AMR_S0 >> t.level[e];
  int64_t p[3];
  for (int d = 0; d < 3; ++d) p[d] = t.origin[3 * (int64_t)e + d] + S / 2;
  const int ax = c_axis[s];
  p[ax] = t.origin[3 * (int64_t)e + ax] + (c_sign[s] > 0 ? S + 1 : -1);
  return d_locate(t, p);
}

__device__ __forceinline__ double shape1d(int order, int i, double xi) {
  if (order == 1) return i == 0 ? __dmul_rn(.5, __dsub_rn(1., xi)) : __dmul_rn(.5, __dadd_rn(1., xi));
  switch (i) {
    case 0: return __dmul_rn(__dmul_rn(.5, xi), __dsub_rn(xi, 1.));
    case 1: return __dmul_rn(__dmul_rn(.5, xi), __dadd_rn(xi, 1.));
    default: return __dmul_rn(__dsub_rn(1., xi), __dadd_rn(1., xi));
  }
}

// QUAD9 / QUAD4 side shape j (fe_lagrange_shape_2D.C node index tables).
__device__ __forceinline__ double side_shape(int ns, int j, double xi, double eta) {
  const int I0[9] = {0, 1, 1, 0, 2, 1, 2, 0, 2}, I1[9] = {0, 0, 1, 1, 0, 2, 1, 2, 2};
  const int order = ns == 9 ? 2 : 1;
  return __dmul_rn(shape1d(order, I0[j], xi), shape1d(order, I1[j], eta));
}

__global__ void k_node_dofs(int64_t n_active, int npe, int n_vars, const int32_t *conn, const int32_t *elem_dofs,
                            int32_t *node_dof) {
  const int64_t total = n_active * npe * n_vars;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = i / (npe * n_vars);
    const int r = (int)(i - a * npe * n_vars), v = r / npe, k = r - v * npe;
    node_dof[(int64_t)conn[a * npe + k] * n_vars + v] = elem_dofs[a * npe * n_vars + v * npe + k];
  }
}

// The visit (v, a, s): whether it applies, and its parent-side data.
struct Visit {
  int32_t e, P;
  int32_t pd[9];
  int64_t L0[3], u[3], w[3], uu, ww;
};

__device__ bool visit(const TreeArgs &t, int64_t i, Visit &x, int &v, int64_t &a, int &s) {
  v = (int)(i / (t.n_active * 6));
  const int64_t r = i - (int64_t)v * t.n_active * 6;
  a = r / 6;
  s = (int)(r - a * 6);
  x.e = t.active[a];
  x.P = t.parent[x.e];
  if (x.P < 0) return false;
  const int c = x.e - t.first_child[x.P];
  bool on = false;
  for (int k = 0; k < 4; ++k) on |= c_hex8[s][k] == c;
  if (!on) return false;  // faces inside the parent meet siblings
  const int32_t nb = d_across(t, x.e, s);
  if (nb < 0 || t.level[nb] >= t.level[x.e]) return false;
  for (int j = 0; j < t.ns; ++j) {
    const int32_t pn = t.tconn[(int64_t)x.P * t.npe + c_sides[s][j]];
    x.pd[j] = t.node_dof[(int64_t)pn * t.n_vars + v];
  }
  const int64_t *L0 = t.node_lat + 3 * (int64_t)t.tconn[(int64_t)x.P * t.npe + c_sides[s][0]];
  const int64_t *L1 = t.node_lat + 3 * (int64_t)t.tconn[(int64_t)x.P * t.npe + c_sides[s][1]];
  const int64_t *L3 = t.node_lat + 3 * (int64_t)t.tconn[(int64_t)x.P * t.npe + c_sides[s][3]];
  x.uu = x.ww = 0;
  for (int d = 0; d < 3; ++d) {
    x.L0[d] = L0[d];
    x.u[d] = L1[d] - L0[d];
    x.w[d] = L3[d] - L0[d];
    x.uu += x.u[d] * x.u[d];
    x.ww += x.w[d] * x.w[d];
  }
  return true;
}

// position of visit (v, a, s) and side node k in libMesh's loop order
__device__ __forceinline__ unsigned long long order_key(const TreeArgs &t, int v, int64_t a, int s, int k) {
  return (((unsigned long long)v * (unsigned long long)t.n_active + (unsigned long long)a) * 6ull + (unsigned)s) *
             16ull + (unsigned)k;
}

template <bool WRITE>
__global__ void k_visits(TreeArgs t) {
  const int64_t total = (int64_t)t.n_vars * t.n_active * 6;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    Visit x;
    int v, s;
    int64_t a;
    if (!visit(t, i, x, v, a, s)) continue;
    for (int k = 0; k < t.ns; ++k) {
      const int32_t my_node = t.tconn[(int64_t)x.e * t.npe + c_sides[s][k]];
      const int32_t my_dof = t.node_dof[(int64_t)my_node * t.n_vars + v];
      bool self = false;
      for (int j = 0; j < t.ns; ++j) self |= x.pd[j] == my_dof;
      if (self) continue;
      if (my_dof < 0 || my_dof >= t.n_dofs) {
        atomicCAS(t.status, 0, (int)LMG_ERR_BOUNDS);
        continue;
      }
      const unsigned long long key = order_key(t, v, a, s, k);
      if (!WRITE) {
        atomicMin(&t.claim[my_dof], key);
        continue;
      }
      if (t.claim[my_dof] != key) continue;
      const int64_t *Lp = t.node_lat + 3 * (int64_t)my_node;
      int64_t pu = 0, pw = 0;
      for (int d = 0; d < 3; ++d) {
        pu += (Lp[d] - x.L0[d]) * x.u[d];
        pw += (Lp[d] - x.L0[d]) * x.w[d];
      }
      const double xi = __dadd_rn(-1., __ddiv_rn(__dmul_rn(2., (double)pu), (double)x.uu));
      const double eta = __dadd_rn(-1., __ddiv_rn(__dmul_rn(2., (double)pw), (double)x.ww));
      // the row's entries in ascending column order (a std::map row), by insertion
      int n = 0;
      int32_t rc[9];
      double rv[9];
      for (int j = 0; j < t.ns; ++j) {
        const double phi = side_shape(t.ns, j, xi, eta);
        if (fabs(phi) > 1.e-5 && fabs(phi) < .999) {
          int q = n++;
          for (; q > 0 && rc[q - 1] > x.pd[j]; --q) {
            rc[q] = rc[q - 1];
            rv[q] = rv[q - 1];
          }
          rc[q] = x.pd[j];
          rv[q] = phi;
        }
      }
      for (int q = 0; q < n; ++q) {
        t.col[(int64_t)my_dof * AMR_ROW_WIDTH + q] = rc[q];
        t.val[(int64_t)my_dof * AMR_ROW_WIDTH + q] = rv[q];
      }
      t.cnt[my_dof] = n;
    }
  }
}

__global__ void k_rows_init(int64_t n, unsigned long long *claim, int32_t *cnt) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    claim[i] = ~0ull;
    cnt[i] = -1;
  }
}

template <typename T>
cudaError_t up(T *&d, const T *h, size_t n) {
  cudaError_t e = cudaMalloc((void **)&d, (n ? n : 1) * sizeof(T));
  if (e == cudaSuccess && n) e = cudaMemcpy(d, h, n * sizeof(T), cudaMemcpyHostToDevice);
  return e;
}

}  // namespace

std::string amr_raw_rows_device(const HostMesh &m, int device, int n_vars, const int32_t *elem_dofs, int64_t n_dofs,
                                std::vector<int32_t> &cnt, std::vector<int32_t> &col, std::vector<double> &val) {
  if (!m.amr.on) {  // no hanging nodes
    cnt.assign((size_t)n_dofs, -1);
    col.clear();
    val.clear();
    return "";
  }
  if (m.elem_type != LMG_HEX8 && m.elem_type != LMG_HEX27) return "device rows: HEX8 or HEX27 meshes";
  if (cudaSetDevice(device) != cudaSuccess) return "device rows: no device";
  const AmrTree &tr = m.amr;
  TreeArgs t{};
  t.nx = tr.nx;
  t.ny = tr.ny;
  t.nz = tr.nz;
  t.npe = m.npe;
  t.n_vars = n_vars;
  t.n_active = (int64_t)tr.active.size();
  t.n_dofs = n_dofs;
  int sides[6][9] = {}, hex8[6][4], vb[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                                {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
  const int axis[6] = {2, 1, 0, 1, 0, 2}, sign[6] = {-1, -1, 1, 1, -1, 1};
  for (int s = 0; s < 6; ++s) {
    t.ns = side_nodes(m.elem_type, s, sides[s]);
    side_nodes(LMG_HEX8, s, hex8[s]);
  }
  const int64_t n_nodes = (int64_t)tr.node_lat.size() / 3;
  int32_t *d_tconn = nullptr, *d_parent = nullptr, *d_fc = nullptr, *d_active = nullptr, *d_conn = nullptr,
          *d_ed = nullptr, *d_nd = nullptr, *d_cnt = nullptr, *d_col = nullptr;
  int8_t *d_level = nullptr;
  int64_t *d_origin = nullptr, *d_lat = nullptr;
  double *d_val = nullptr;
  unsigned long long *d_claim = nullptr;
  int *d_status = nullptr;
  std::string err;
  cudaError_t e = cudaSuccess;
  auto ok = [&](cudaError_t x) {
    if (e == cudaSuccess) e = x;
    return e == cudaSuccess;
  };
  const int64_t nl = (int64_t)m.npe * n_vars;
  if (ok(cudaMemcpyToSymbol(c_sides, sides, sizeof(sides))) && ok(cudaMemcpyToSymbol(c_hex8, hex8, sizeof(hex8))) &&
      ok(cudaMemcpyToSymbol(c_vbits, vb, sizeof(vb))) && ok(cudaMemcpyToSymbol(c_axis, axis, sizeof(axis))) &&
      ok(cudaMemcpyToSymbol(c_sign, sign, sizeof(sign))) && ok(up(d_tconn, tr.conn.data(), tr.conn.size())) &&
      ok(up(d_parent, tr.parent.data(), tr.parent.size())) &&
      ok(up(d_fc, tr.first_child.data(), tr.first_child.size())) &&
      ok(up(d_level, tr.level.data(), tr.level.size())) && ok(up(d_origin, tr.origin.data(), tr.origin.size())) &&
      ok(up(d_lat, tr.node_lat.data(), tr.node_lat.size())) &&
      ok(up(d_active, tr.active.data(), tr.active.size())) && ok(up(d_conn, m.conn.data(), m.conn.size())) &&
      ok(up(d_ed, elem_dofs, (size_t)(t.n_active * nl))) &&
      ok(cudaMalloc((void **)&d_nd, sizeof(int32_t) * (size_t)(n_nodes * n_vars))) &&
      ok(cudaMemset(d_nd, 0xff, sizeof(int32_t) * (size_t)(n_nodes * n_vars))) &&
      ok(cudaMalloc((void **)&d_claim, sizeof(unsigned long long) * (size_t)n_dofs)) &&
      ok(cudaMalloc((void **)&d_cnt, sizeof(int32_t) * (size_t)n_dofs)) &&
      ok(cudaMalloc((void **)&d_col, sizeof(int32_t) * (size_t)n_dofs * AMR_ROW_WIDTH)) &&
      ok(cudaMalloc((void **)&d_val, sizeof(double) * (size_t)n_dofs * AMR_ROW_WIDTH)) &&
      ok(cudaMalloc((void **)&d_status, sizeof(int))) && ok(cudaMemset(d_status, 0, sizeof(int)))) {
    t.tconn = d_tconn;
    t.parent = d_parent;
    t.first_child = d_fc;
    t.level = d_level;
    t.origin = d_origin;
    t.node_lat = d_lat;
    t.active = d_active;
    t.node_dof = d_nd;
    t.claim = d_claim;
    t.cnt = d_cnt;
    t.col = d_col;
    t.val = d_val;
    t.status = d_status;
    const int threads = 256;
    auto blocks = [&](int64_t n) { return (int)std::min<int64_t>((n + threads - 1) / threads, 65536); };
    k_node_dofs<<<blocks(t.n_active * nl), threads>>>(t.n_active, m.npe, n_vars, d_conn, d_ed, d_nd);
    k_rows_init<<<blocks(n_dofs), threads>>>(n_dofs, d_claim, d_cnt);
    const int64_t visits = (int64_t)n_vars * t.n_active * 6;
    k_visits<false><<<blocks(visits), threads>>>(t);
    k_visits<true><<<blocks(visits), threads>>>(t);
    int status = 0;
    if (ok(cudaGetLastError()) && ok(cudaDeviceSynchronize()) &&
        ok(cudaMemcpy(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost))) {
      if (status) {
        err = "constraints: dof out of range";
      } else {
        cnt.resize((size_t)n_dofs);
        col.resize((size_t)n_dofs * AMR_ROW_WIDTH);
        val.resize((size_t)n_dofs * AMR_ROW_WIDTH);
        ok(cudaMemcpy(cnt.data(), d_cnt, sizeof(int32_t) * cnt.size(), cudaMemcpyDeviceToHost));
        ok(cudaMemcpy(col.data(), d_col, sizeof(int32_t) * col.size(), cudaMemcpyDeviceToHost));
        ok(cudaMemcpy(val.data(), d_val, sizeof(double) * val.size(), cudaMemcpyDeviceToHost));
      }
    }
  }
  if (e != cudaSuccess && err.empty()) err = std::string("device rows: ") + cudaGetErrorString(e);
  for (void *p : {(void *)d_tconn, (void *)d_parent, (void *)d_fc, (void *)d_active, (void *)d_conn, (void *)d_ed,
                  (void *)d_nd, (void *)d_cnt, (void *)d_col, (void *)d_level, (void *)d_origin, (void *)d_lat,
                  (void *)d_val, (void *)d_claim, (void *)d_status})
    if (p) cudaFree(p);
  return err;
}

}  // namespace lmg
