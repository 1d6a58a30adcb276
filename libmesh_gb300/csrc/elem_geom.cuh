// Element geometry shared by the element kernels (elements.cu, tc.cu): the
// FP64 map of compute_affine_map / compute_single_point_map, the Lame
// constants of the elasticity form and the FP64 load-vector contribution of
// one quadrature point.  One definition, so that every kernel using them gets
// the same bits.
#pragma once

#include <cuda_runtime.h>

namespace lmg {

// Jacobian at one point from the mapping shape derivatives gd [n_geo][3] and
// element coordinates X [n_geo][3]; returns detJ and G[m][d] = dxi_m / dx_d.
__device__ __forceinline__ double invert_map(const double J[9], double G[9]);

__device__ __forceinline__ double jacobian(const double *X, const double *gd, int n_geo,
                                           double G[9]) {
  double J[9];  // J[m*3+d] = d x_d / d xi_m
#pragma unroll
  for (int i = 0; i < 9; ++i) J[i] = 0.0;
  for (int a = 0; a < n_geo; ++a) {
    const double x = X[3 * a], y = X[3 * a + 1], z = X[3 * a + 2];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const double g = gd[3 * a + m];
      J[3 * m + 0] += x * g;
      J[3 * m + 1] += y * g;
      J[3 * m + 2] += z * g;
    }
  }
  return invert_map(J, G);
}

// The constant map of an affine element (compute_affine_map's value) from the
// edge vectors of its vertices: tets v1 - v0, v2 - v0, v3 - v0; hexahedra
// (v1 - v0) / 2, (v3 - v0) / 2, (v4 - v0) / 2 (reference edge length 2);
// prisms v1 - v0, v2 - v0, (v3 - v0) / 2.  N, the element's node count,
// identifies the type (4, 10 tets; 8, 27 hexahedra; 6 prisms).
template <int N>
__device__ __forceinline__ double jacobian_affine(const double *X, double G[9]) {
  constexpr bool hex = (N == 8 || N == 27);
  constexpr int v[3] = {1, hex ? 3 : 2, hex ? 4 : 3};
  constexpr double sc[3] = {hex ? 0.5 : 1.0, hex ? 0.5 : 1.0, (hex || N == 6) ? 0.5 : 1.0};
  double J[9];
#pragma unroll
  for (int m = 0; m < 3; ++m)
#pragma unroll
    for (int d = 0; d < 3; ++d) J[3 * m + d] = sc[m] * (X[3 * v[m] + d] - X[d]);
  return invert_map(J, G);
}

__device__ __forceinline__ double invert_map(const double J[9], double G[9]) {
  const double xxi = J[0], yxi = J[1], zxi = J[2];
  const double xet = J[3], yet = J[4], zet = J[5];
  const double xze = J[6], yze = J[7], zze = J[8];
  const double c0 = yet * zze - zet * yze, c1 = zet * xze - xet * zze, c2 = xet * yze - yet * xze;
  const double det = xxi * c0 + yxi * c1 + zxi * c2;
  const double inv = 1.0 / det;
  G[0] = c0 * inv;
  G[1] = c1 * inv;
  G[2] = c2 * inv;
  G[3] = (zxi * yze - yxi * zze) * inv;
  G[4] = (xxi * zze - zxi * xze) * inv;
  G[5] = (yxi * xze - xxi * yze) * inv;
  G[6] = (yxi * zet - zxi * yet) * inv;
  G[7] = (zxi * xet - xxi * zet) * inv;
  G[8] = (xxi * yet - yxi * xet) * inv;
  return det;
}

// Lamé constants of libMesh's elasticity_tensor with Young's modulus E.
__device__ __forceinline__ void lame(double E, double nu, double &lam, double &mu) {
  lam = (E * nu) / ((1. + nu) * (1. - 2. * nu));
  mu = E / (2. * (1. + nu));
}

// Load vector of one element, F_a^v = sum_q (JxW_q f^v(x_q)) phi_a(q) with
// f^v(x_q) = sum_b phi_b(q) f_b^v (the FE interpolation of the nodal load),
// both sums in order with explicit fused multiply-adds, by one warp: first
// lane (q, v) forms f^v(x_q) into fq [Q][NV], then lane (a, v) the sum over q.
// ph = phi [Q][N], f = nodal load [N][NV], jxw [Q] (stride jstride), fq scratch
// [Q][NV]; out(a, v, value) receives each entry.
template <int N, int NV, typename Out>
__device__ __forceinline__ void element_load(const double *ph, const double *f, const double *jxw, int jstride, int Q,
                                             double *fq, int lane, Out &&out) {
  for (int idx = lane; idx < Q * NV; idx += 32) {
    const int q = idx / NV, v = idx - q * NV;
    double s = 0.0;
    for (int b = 0; b < N; ++b) s = fma(ph[q * N + b], f[b * NV + v], s);
    fq[idx] = s;
  }
  __syncwarp();
  for (int idx = lane; idx < N * NV; idx += 32) {
    const int a = idx / NV, v = idx - a * NV;
    double acc = 0.0;
    for (int q = 0; q < Q; ++q) acc = fma(jxw[q * jstride] * fq[q * NV + v], ph[q * N + a], acc);
    out(a, v, acc);
  }
  __syncwarp();
}

}  // namespace lmg
